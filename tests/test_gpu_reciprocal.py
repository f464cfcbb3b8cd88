"""The device reciprocal of the flux kernels (rcp.approx.ftz.f64 estimate refined by two Newton-Raphson steps,
sdg_device.cuh `rcp`) against IEEE 1/x: within 1 ulp wherever x and 1/x are normal doubles, over the whole
exponent range and at the densities and pressures a flow has."""
import ctypes

import numpy as np
import pytest

from subrosadg_gb300 import _abi

pytestmark = pytest.mark.gpu


def _device_reciprocal(x):
    lib = _abi.load()
    x = np.ascontiguousarray(x, np.float64)
    out = np.empty_like(x)
    p = ctypes.POINTER(ctypes.c_double)
    _abi.check(lib.sdg_probe_reciprocal(0, x.ctypes.data_as(p), out.ctypes.data_as(p), x.size))
    return out


def _ulps(a, b):
    """Distance in units in the last place between doubles of the same sign."""
    ia, ib = a.view(np.int64), b.view(np.int64)
    return np.abs(ia - ib)


def test_reciprocal_within_one_ulp_over_the_normal_range():
    rng = np.random.default_rng(17)
    exps = rng.integers(-1021, 1022, 200_000)
    mant = rng.uniform(1.0, 2.0, exps.size)
    x = np.ldexp(mant, exps)
    x = np.concatenate([x, -x[:1000], np.ldexp(1.0, np.arange(-1021, 1022)),      # powers of two: exact
                        np.nextafter(1.0, [0.0, 2.0]), rng.uniform(1e-3, 1e3, 50_000)])  # near 1, flow values
    r = _device_reciprocal(x)
    ref = 1.0 / x
    assert np.all(np.isfinite(r))
    assert np.all(np.sign(r) == np.sign(ref))
    err = _ulps(np.abs(r), np.abs(ref))
    assert err.max() <= 1, f"max {err.max()} ulp at x = {x[np.argmax(err)]!r}"
    exact = np.ldexp(1.0, -np.arange(-1021, 1022))
    np.testing.assert_array_equal(r[201_000:201_000 + exact.size], exact)


def test_reciprocal_rejects_bad_arguments():
    lib = _abi.load()
    p = ctypes.POINTER(ctypes.c_double)
    x = np.ones(4)
    assert lib.sdg_probe_reciprocal(0, x.ctypes.data_as(p), x.ctypes.data_as(p), 0) == _abi.SDG_ERR_INVALID_ARGUMENT
    assert lib.sdg_probe_reciprocal(0, None, x.ctypes.data_as(p), 4) == _abi.SDG_ERR_INVALID_ARGUMENT
