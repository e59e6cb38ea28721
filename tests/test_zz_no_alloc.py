"""icm_gpu_equity_noalloc: the entry point for callers that cannot allocate
device memory (hosts that forbid device allocation after start-up, processes
whose device memory belongs to another allocator's pool).  Its device
data lives in the library's static scratch array, so each call overwrites
the last; two calls in a row must both agree with icm_equity.

This file runs last (pytest collects it after the other test files) so that
a failure here cannot hide another test's result in a run that stops at the
first failure.  It passes alone in a fresh process and after the others."""
import ctypes

import numpy as np
import pytest

from tests.conftest import max_rel
from icm_gb300 import workloads as W

pytestmark = pytest.mark.gpu

_dp = ctypes.POINTER(ctypes.c_double)


def _noalloc(L, S, P, Q=256):
    S = np.ascontiguousarray(S, dtype=np.float64)
    P = np.ascontiguousarray(P, dtype=np.float64)
    out = np.full(len(S), np.nan)
    rc = L.icm_gpu_equity_noalloc(len(S), S.ctypes.data_as(_dp), Q, P.ctypes.data_as(_dp), len(P),
                                  out.ctypes.data_as(_dp))
    return rc, out


@pytest.mark.parametrize("case", ["plain_small", "dropin_4096", "truncated_3000", "tiny"])
def test_noalloc_matches_icm_equity_on_two_calls(gpu_icm, case):
    from icm_gb300._lib import lib
    L = lib()
    if case == "plain_small":
        S, P = W.plain_small()
    elif case == "dropin_4096":
        S, P, _ = W.dropin(n=4096)
    elif case == "truncated_3000":   # k < n: truncated (coefficient-FFT) levels above the crossover
        rng = np.random.default_rng(30)
        S, P = 1e4 * np.exp(rng.standard_normal(3000)), W.geometric_payout(450, 0.99)
    else:
        S, P = np.array([3.0, 1.0, 2.0]), np.array([0.7, 0.3])
    ref = gpu_icm.equity(S, P)
    for _ in range(2):    # the second call reuses scratch the first one filled
        rc, out = _noalloc(L, S, P)
        assert rc == 0, L.icm_gpu_last_error().decode()
        assert max_rel(out, ref) < 1e-12


def test_noalloc_rejects_sizes_beyond_its_limit(gpu_icm):
    from icm_gb300._lib import lib
    L = lib()
    S = np.linspace(1.0, 2.0, 4097)
    rc, out = _noalloc(L, S, np.array([1.0]))
    assert rc == -1
    assert "4096" in L.icm_gpu_last_error().decode()
    rc, out = _noalloc(L, S[:100], np.array([1.0]), Q=5000)
    assert rc == -1
    assert "limit" in L.icm_gpu_last_error().decode()
