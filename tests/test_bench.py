"""bench.py's host-side arithmetic: the reference's canonical work per solve
(restated from its tree geometry and FFT-tier counts) for the measured
configurations, against the figures the reference's cost model gives for
them: drop-in 8.93e10 flop / 1.36e10 B, n = k = 2^20 2.25e12 / 3.24e11,
n = 2^20, k = 1000 6.46e11 / 8.5e10, n = 16384, k = 2000 1.22e10 / 2.0e9."""
import pytest

import bench


@pytest.mark.parametrize("n,k,W,D", [(65536, 65536, 8.93e10, 1.36e10), (1 << 20, 1 << 20, 2.25e12, 3.24e11),
                                     (1 << 20, 1000, 6.46e11, 8.5e10), (16384, 2000, 1.22e10, 2.0e9)])
def test_canonical_work(n, k, W, D):
    w, d = bench.canonical_work(n, k, bench.REF_B[(n, k)])
    assert abs(w / W - 1) < 0.005 and abs(d / D - 1) < 0.011


def test_canonical_rates():
    r = bench.canonical_rates(65536, 65536, 20.0, 1.25)
    assert r["B_ref"] == 64 and r["achieved_fp64"] == pytest.approx(8.931e10 / (0.02 * 1.25e12), rel=1e-3)
    assert bench.canonical_rates(1000, 10, 1.0, 1.25) is None
