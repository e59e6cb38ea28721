"""Seeded synthetic tournaments for parity tests and benchmarks.

Every generator is driven by splitmix64 (the generator the reference uses for
its golden vectors, ``web/verify/gen_reference.c:19-32``) in numpy uint64
arithmetic, so the same seed gives the same stacks on x86 and Arm hosts.
Normal deviates use Box-Muller; Gamma(2, theta) is the sum of two
exponentials.  Shapes follow the five workloads the reference's scope lists:

* ``plain_small``   n=1024, k=100, integer stacks U[1,10000], linear payouts
* ``dropin``        n=k=65536, log-uniform stacks over [1,1e9], quadratic payouts,
                    plus 64 distinct subset targets
* ``gpu_scale``     n=1,048,576, stacks 1e4*lognormal(0,1.5); k=n linear or
                    k=1000 geometric (0.97)
* ``batched``       4096 tournaments, n log-uniform in [9,20000],
                    k=min(n,ceil(0.15 n)), stacks 1e4*lognormal(0,1),
                    geometric payouts (0.8)
* ``vjp``           n=16384, k=2000, stacks Gamma(2,5000), linear/quadratic payouts
* ``b200_heatmap``  the inputs of the reference's published B200 timings:
                    stacks 1 + 99 U(0,1), unnormalised payout n - m

All payouts are normalised to sum 1 unless stated otherwise.
"""
from __future__ import annotations

import math

import numpy as np

_GAMMA = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)
SEED = 0x1CEB00DA


class SplitMix64:
    """splitmix64 stream; ``uniform`` matches gen_reference.c's ``uni``."""

    def __init__(self, seed: int = SEED):
        self.state = np.uint64(seed)

    def next_u64(self, count: int) -> np.ndarray:
        with np.errstate(over="ignore"):
            steps = np.arange(1, count + 1, dtype=np.uint64)
            z = self.state + steps * _GAMMA
            self.state = self.state + np.uint64(count) * _GAMMA
            z = (z ^ (z >> np.uint64(30))) * _M1
            z = (z ^ (z >> np.uint64(27))) * _M2
            return z ^ (z >> np.uint64(31))

    def uniform(self, count: int, lo: float = 0.0, hi: float = 1.0) -> np.ndarray:
        u = (self.next_u64(count) >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)
        return lo + u * (hi - lo)

    def integers(self, count: int, lo: int, hi: int) -> np.ndarray:
        """Uniform integers in [lo, hi] (inclusive)."""
        u = self.uniform(count)
        return lo + np.floor(u * (hi - lo + 1)).astype(np.int64)

    def normal(self, count: int) -> np.ndarray:
        u1 = 1.0 - self.uniform(count)          # (0, 1]
        u2 = self.uniform(count)
        return np.sqrt(-2.0 * np.log(u1)) * np.cos(2.0 * math.pi * u2)

    def exponential(self, count: int) -> np.ndarray:
        return -np.log(1.0 - self.uniform(count))


def normalise(p: np.ndarray) -> np.ndarray:
    return p / p.sum()


def linear_payout(k: int) -> np.ndarray:
    return normalise(np.arange(k, 0, -1, dtype=np.float64))


def quadratic_payout(k: int) -> np.ndarray:
    return normalise(np.arange(k, 0, -1, dtype=np.float64) ** 2)


def geometric_payout(k: int, ratio: float) -> np.ndarray:
    return normalise(ratio ** np.arange(k, dtype=np.float64))


def plain_small(n: int = 1024, k: int = 100, seed: int = SEED):
    rng = SplitMix64(seed)
    S = rng.integers(n, 1, 10000).astype(np.float64)
    return S, linear_payout(k)


def dropin(n: int = 65536, k: int | None = None, n_targets: int = 64, seed: int = SEED + 2):
    k = n if k is None else k
    rng = SplitMix64(seed)
    S = 10.0 ** rng.uniform(n, 0.0, 9.0)
    # distinct targets: partial Fisher-Yates driven by the same stream
    idx = np.arange(n)
    r = rng.uniform(n_targets)
    for t in range(n_targets):
        j = t + int(r[t] * (n - t))
        idx[t], idx[j] = idx[j], idx[t]
    targets = np.sort(idx[:n_targets]).astype(np.int32)
    return S, quadratic_payout(k), targets


def gpu_scale(n: int = 1 << 20, shape: str = "linear", seed: int = SEED + 3):
    rng = SplitMix64(seed)
    S = 1e4 * np.exp(1.5 * rng.normal(n))
    if shape == "linear":
        return S, linear_payout(n)
    return S, geometric_payout(min(1000, n), 0.97)


def batched(count: int = 4096, n_lo: int = 9, n_hi: int = 20000, seed: int = SEED + 4):
    """List of (stacks, payout) for independent tournaments."""
    rng = SplitMix64(seed)
    ns = np.rint(np.exp(rng.uniform(count, math.log(n_lo), math.log(n_hi)))).astype(np.int64)
    out = []
    for n in ns:
        n = int(n)
        k = min(n, int(math.ceil(0.15 * n)))
        S = 1e4 * np.exp(rng.normal(n))
        out.append((S, geometric_payout(k, 0.8)))
    return out


def vjp(n: int = 16384, k: int = 2000, payout: str = "linear", seed: int = SEED + 5):
    rng = SplitMix64(seed)
    S = 5000.0 * (rng.exponential(n) + rng.exponential(n))
    P = linear_payout(k) if payout == "linear" else quadratic_payout(k)
    cot = rng.normal(n)
    return S, P, cot


def b200_heatmap(n: int = 65536, k: int | None = None, seed: int = SEED + 6):
    """The inputs of the reference's published B200 timings
    (tools/heatmap_gpu.cu:15-25): stacks 1 + 99 U(0,1), payout n - m
    (unnormalised), m < k.  The reference draws U from the C library's rand()
    seeded with 42 + n; here it is splitmix64 (same distribution; the tree's
    work depends on the stacks only through their spread)."""
    k = n if k is None else k
    rng = SplitMix64(seed)
    S = 1.0 + 99.0 * rng.uniform(n)
    return S, (n - np.arange(k)).astype(np.float64)
