"""Inputs of the reference's golden vectors (web/verify/reference.json).

The reference's generator (web/verify/gen_reference.c:19-137) draws every
case from one splitmix64 stream seeded with 0x1CEB00DA, in a fixed case order.
This module restates that generator so tests can rebuild each case's stacks
and payouts exactly; tests/golden/web_reference.json stores only the
reference's equities.  make_golden.py checks the rebuilt stacks against
reference.json bit for bit before writing the fixture.
"""
from __future__ import annotations

import numpy as np

from fractions import Fraction

from icm_gb300.workloads import SplitMix64


def _uni(rng: SplitMix64, count: int, lo: float, hi: float) -> np.ndarray:
    """gen_reference.c's uni(): lo + u*(hi-lo).  The golden file was made by
    a compiler that contracts this into one fused multiply-add, so the sum is
    rounded once, from the exact value."""
    u = rng.uniform(count)
    span = Fraction(hi - lo)
    return np.array([float(Fraction(lo) + Fraction(float(x)) * span) for x in u])

# (name, n, k, Q, kind, pool): gen_reference.c:121-136
CASES = [
    ("headsup", 2, 1, 256, "uniform", 1.0),
    ("ft9", 9, 3, 256, "uniform", 1.0),
    ("sng10", 10, 10, 256, "uniform", 1.0),
    ("mtt45", 45, 7, 256, "loguniform", 45000.0),
    ("mtt200", 200, 27, 512, "loguniform", 200000.0),
    ("mtt1000", 1000, 150, 1024, "loguniform", 1e6),
    ("mtt3000", 3000, 450, 1024, "loguniform", 3e6),
    ("mtt10000", 10000, 1500, 2048, "loguniform", 1e7),
    ("allpaid2000", 2000, 2000, 256, "uniform", 1.0),
    ("ratio1e9", 9, 3, 256, "ratio1e9", 1.0),
    ("ratio1e9_100", 100, 15, 512, "ratio1e9", 1.0),
    ("equal100", 100, 15, 256, "equal", 1.0),
    ("cash6", 6, 2, 256, "uniform", 2000.0),
    ("k1_500", 500, 1, 256, "loguniform", 1.0),
    ("allpaid300", 300, 300, 256, "loguniform", 1.0),
    ("linear27", 27, 5, 256, "uniform", 1.0),
]


def _stacks(rng: SplitMix64, n: int, kind: str) -> np.ndarray:
    if kind == "uniform":
        return _uni(rng, n, 500.0, 200000.0)
    if kind == "equal":
        return np.full(n, 10000.0)
    if kind == "ratio1e9":
        S = np.empty(n)
        S[0], S[1] = 1.0, 1e9
        S[2:] = _uni(rng, n - 2, 1.0, 1e9)
        return S
    # loguniform: per player e = uni(0,6) then uni(1,10) * 10^floor(e),
    # the power built by repeated multiplication as the C code does
    S = np.empty(n)
    for i in range(n):
        e = _uni(rng, 1, 0.0, 6.0)[0]
        m = 1.0
        for _ in range(int(e)):
            m *= 10.0
        S[i] = _uni(rng, 1, 1.0, 10.0)[0] * m
    return S


def _payouts(k: int, pool: float) -> np.ndarray:
    p = 1.0 / (1.0 + 0.5 * np.arange(k, dtype=np.float64))
    s = 0.0
    for v in p:           # sequential sum, as the C loop
        s += v
    return p * (pool / s)


def all_cases():
    """Yield (name, n, k, Q, stacks, payouts) in the reference's order."""
    rng = SplitMix64(0x1CEB00DA)
    for name, n, k, Q, kind, pool in CASES:
        yield name, n, k, Q, _stacks(rng, n, kind), _payouts(k, pool)
