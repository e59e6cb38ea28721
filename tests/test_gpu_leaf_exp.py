"""The leaves' exponential (a table-driven exp on [-700, 0]) against the
host's exp: within one unit in the last place everywhere, 0 below -700
(reference src/cpu/icm.c:2575-2581, the leaf factor's cut-off)."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

_dp = ctypes.POINTER(ctypes.c_double)


def _leaf(gpu_icm, x):
    from icm_gb300._lib import lib
    x = np.ascontiguousarray(x, dtype=np.float64)
    out = np.full(len(x), np.nan)
    assert lib().icm_gb300_leaf_factors(len(x), x.ctypes.data_as(_dp), out.ctypes.data_as(_dp)) == 0
    return out


def _ulps(a, b):
    return np.abs(a.view(np.int64) - b.view(np.int64))


def test_leaf_exp_within_one_ulp(gpu_icm):
    rng = np.random.default_rng(11)
    ln2_128 = np.log(2.0) / 128
    x = np.concatenate([
        -700.0 * rng.random(1 << 20),                       # the whole domain
        -rng.random(1 << 16) * 1e-3,                        # near 0
        -np.logspace(-300, 0, 4096),                        # tiny arguments
        -700.0 + rng.random(4096) * 1e-3,                   # near the cut-off
        -np.arange(1, 700 * 128) * ln2_128,                 # reduction boundaries
        -(np.arange(1, 4096) + 0.5) * ln2_128,              # the largest |r|
        [0.0, -0.0, -700.0, -1e-300, -5e-324],
    ])
    got = _leaf(gpu_icm, x)
    ref = np.exp(x)
    u = _ulps(got, ref)
    assert u.max() <= 1, (u.max(), x[np.argmax(u)])
    assert np.mean(u == 0) > 0.9
    assert got[-5] == 1.0 and got[-4] == 1.0


def test_leaf_exp_cut_off(gpu_icm):
    x = np.array([-700.0000001, -701.0, -745.0, -1e6, -np.inf])
    assert np.all(_leaf(gpu_icm, x) == 0.0)
